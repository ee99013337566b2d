set output "hist_sp_MOTIF00003.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-52.2817:18.834]
set yrange [0:7775]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00003.dat" using 1:2 title 'MOTIF00003 (sp)' with boxes
