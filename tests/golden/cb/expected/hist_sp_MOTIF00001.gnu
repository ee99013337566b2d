set output "hist_sp_MOTIF00001.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-61.1576:22.3747]
set yrange [0:8637]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00001.dat" using 1:2 title 'MOTIF00001 (sp)' with boxes
