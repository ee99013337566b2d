set output "hist_sp_MOTIF00005.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-58.8019:18.7062]
set yrange [0:7658]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00005.dat" using 1:2 title 'MOTIF00005 (sp)' with boxes
