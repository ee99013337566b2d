set output "hist_sp_MOTIF00000.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-52.4869:17.989]
set yrange [0:7194]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00000.dat" using 1:2 title 'MOTIF00000 (sp)' with boxes
